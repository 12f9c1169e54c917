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


@pytest.mark.parametrize("n", [231, 232, 233])
def test_eigen_solve_tridiagonal_limit(ctx, n):
    """Up to 232 the eigen-solve runs Householder + bisection + inverse
    iteration; from 233 the Jacobi solver.  Both against LAPACK."""
    a = np.random.default_rng(1000 + n).standard_normal((n, n))
    a = a + a.T
    w, v = ctx.eigen_solve(a)
    wr = np.linalg.eigvalsh(a)
    sc = np.abs(wr).max()
    np.testing.assert_allclose(w, wr, rtol=0, atol=1e-12 * sc)
    assert np.max(np.abs(a @ v - v * w)) < 1e-11 * sc
    assert np.max(np.abs(v.T @ v - np.eye(n))) < 1e-12


def _clustered(n_cl, rng):
    lam = np.concatenate([np.full(10, -3.0) + 1e-12 * np.arange(10), np.linspace(0.0, 1.0, n_cl),
                          5.0 + 1e-9 * np.arange(10), np.repeat([7.0, 8.0], 5)])
    q, _ = np.linalg.qr(rng.standard_normal((lam.size, lam.size)))
    return q @ np.diag(lam) @ q.T, lam


def test_eigen_solve_clustered_and_repeated(ctx):
    """Eigenvalues 1e-12 and 1e-9 apart and exactly repeated ones in a dense
    matrix: orthonormal eigenvectors with small residuals."""
    a, lam = _clustered(100, np.random.default_rng(5))
    w, v = ctx.eigen_solve(a)
    np.testing.assert_allclose(w, np.sort(lam), rtol=0, atol=1e-13 * 8)
    assert np.max(np.abs(a @ v - v * w)) < 1e-13 * 8
    assert np.max(np.abs(v.T @ v - np.eye(lam.size))) < 1e-13


def test_eigen_solve_scf_fock_both_solvers():
    """The orthogonal-basis Fock matrix of (H2O)4/STO-3G at convergence (near-
    degenerate O 1s levels 1e-3 apart): tridiagonal solver and Jacobi agree."""
    import os
    fb = B.flatten(M.cluster_atoms("batch256", "sto-3g", index=20))
    ob = O.OracleBasis(fb)
    r = O.scf(fb, O.SCFOptions.baseline(guess="sad"))
    x = O.symm_ortho(O.tri_to_square(ob.overlap(False)))
    fp = x.T @ O.tri_to_square(r.fock) @ x
    with _lib.Context(0) as c:
        w, v = c.eigen_solve(fp)
    old = os.environ.get("GBHF_EIGEN")
    os.environ["GBHF_EIGEN"] = "jacobi"
    try:
        with _lib.Context(0) as c:
            wj, vj = c.eigen_solve(fp)
    finally:
        if old is None:
            del os.environ["GBHF_EIGEN"]
        else:
            os.environ["GBHF_EIGEN"] = old
    wr = np.linalg.eigvalsh(fp)
    np.testing.assert_allclose(w, wr, rtol=0, atol=1e-12 * 21)
    np.testing.assert_allclose(wj, wr, rtol=0, atol=1e-12 * 21)
    assert np.max(np.abs(np.abs(np.sum(v * vj, axis=0)) - 1.0)) < 1e-9
    assert np.max(np.abs(v.T @ v - np.eye(fp.shape[0]))) < 1e-13


@pytest.mark.parametrize("n", [16, 17, 100, 232])
def test_tridiagonalisation_cluster_and_single_cta(ctx, n):
    """The 8-CTA cluster tridiagonalisation (the default) and the one-CTA form
    (GBHF_EIGEN=single-cta) both give LAPACK's spectrum and orthonormal vectors."""
    import os
    a = np.random.default_rng(2000 + n).standard_normal((n, n))
    a = a + a.T
    wr = np.linalg.eigvalsh(a)
    sc = np.abs(wr).max()
    w, v = ctx.eigen_solve(a)
    old = os.environ.get("GBHF_EIGEN")
    os.environ["GBHF_EIGEN"] = "single-cta"
    try:
        with _lib.Context(0) as c:
            w1, v1 = c.eigen_solve(a)
    finally:
        if old is None:
            del os.environ["GBHF_EIGEN"]
        else:
            os.environ["GBHF_EIGEN"] = old
    for ww, vv in ((w, v), (w1, v1)):
        np.testing.assert_allclose(ww, wr, rtol=0, atol=1e-12 * sc)
        assert np.max(np.abs(a @ vv - vv * ww)) < 1e-11 * sc
        assert np.max(np.abs(vv.T @ vv - np.eye(n))) < 1e-12
