"""Pin the oracle against the known-answer data the reference carries.

* Boys function: the Mamedov (2004) table quoted in
  Science/QuantumChemistry/NumericalTools/Boys.hs:27-39 ("Eq(3)" column; the
  m=20, x=30 entry is printed there as 1.37585444267909e-3, a misprint of
  e-13: F_20(30) ~ 39!!/(2^21) sqrt(pi/30^41) ~ 1.4e-13, and the reference's
  own "ours" column in the same comment reads 1.3758e-13).
* Gauss elimination: the system q1/v1 of
  NumericalTools/GaussElimination.hs:115-119, solution (1, -2, 3).
* 256-point Gauss-Legendre table of PointsWeights.hs: hash + deviation
  recorded in tests/golden/quadrature256.json (made by make_golden.py).
* Textbook energies of the STO-3G systems the reference's driver follows
  (Szabo & Ostlund, cited in HartreeFock/HartreeFock.hs:20-21).
"""
import hashlib
import re

import numpy as np
import pytest

import oracle as O
from conftest import REFERENCE, golden
from gbhf import basis as B

MAMEDOV = [(8, 16, 4.02308592502660e-07), (15, 27, 1.08359515555596e-11), (20, 30, 1.37585444267909e-13),
           (25, 13, 8.45734447905704e-08), (31, 34, 2.90561943091301e-16), (11, 38, 4.04561442253925e-12),
           (42, 32, 5.02183610419087e-16), (75, 30, 1.01429517438537e-15), (100, 33, 3.42689684943483e-17),
           (20, 1.4e-3, 2.43577075309547e-02), (45, 6.4e-5, 1.09883228385254e-02),
           (100, 2.6e-7, 4.97512309732144e-03)]


@pytest.mark.parametrize("m,x,v", MAMEDOV)
def test_boys_exact_matches_mamedov_table(m, x, v):
    assert O.boys_exact(m, x) == pytest.approx(v, rel=1e-13)


@pytest.mark.parametrize("m,x,v", MAMEDOV)
def test_boys_reference_quadrature_matches_mamedov_table(m, x, v):
    # the reference's own boysF (Kummer integral, 256-point rule)
    assert O.boys_ref(m, x) == pytest.approx(v, rel=1e-13)


def test_reference_grid_error_bounds():
    """generateGridBoys 0.1 versus the exact function: F_0 exact, F_1 carries the
    quadrature error of the t^(1/2) integrand (<= 3.1e-9 absolute), m >= 2 below 1e-13."""
    g = O.boys_ref_grid()
    xs = np.arange(1001) * 0.1
    for m in range(15):
        ex = np.array([O.boys_exact(m, x) for x in xs[::7]])
        err = np.max(np.abs(g[m, ::7] - ex))
        bound = {0: 1e-15, 1: 3.1e-9, 2: 4e-14}.get(m, 1e-15)
        assert err <= bound, (m, err)


def test_gauss_elimination_known_answer():
    x = O.gauss_elem([[4.0, -2.0, 1.0], [-2.0, 4.0, -2.0], [1.0, -2.0, 4.0]], [11.0, -16.0, 17.0])
    np.testing.assert_allclose(x, [1.0, -2.0, 3.0], rtol=0, atol=1e-14)


def test_gauss_elimination_failure_rules():
    # a row without any |entry| > 1e-6 after elimination -> Nothing
    assert O.gauss_elem([[1.0, 2.0], [2.0, 4.0]], [1.0, 2.0]) is None
    assert O.gauss_elem([[np.nan, 0.0], [0.0, 1.0]], [1.0, 1.0]) is None
    assert O.gauss_elem([[0.0, 1.0], [1.0, 0.0]], [1.0, 1.0]) is None   # zero pivot -> Inf


def _pw_table():
    src = (REFERENCE / "Science/QuantumChemistry/NumericalTools/PointsWeights.hs").read_text()

    def get(name):
        m = re.search(name + r" = U.fromList \[([^\]]*)\]", src)
        return np.array([float(v) for v in m.group(1).split(",")])
    return get("points256"), get("weights256")


def test_gauss_legendre_nodes_match_reference_table():
    fix = golden("quadrature256.json")
    x, w = O.gauss_legendre(256)
    assert x.size == fix["n_positive_nodes"] == 128
    # Gauss-Legendre exactness: integrate x^k on [-1,1] for k < 2n
    for k in (0, 2, 10, 100, 254):
        assert 2 * np.sum(w * x ** k) == pytest.approx(2.0 / (k + 1), rel=1e-13)
    if REFERENCE is not None and (REFERENCE / "Science").exists():
        px, pw = _pw_table()
        h = hashlib.sha256(np.asarray(px, ">f8").tobytes() + np.asarray(pw, ">f8").tobytes()).hexdigest()
        assert h == fix["reference_sha256"]
        assert np.max(np.abs(x - px)) == 0.0
        assert np.max(np.abs(w - pw)) <= 4e-18
    else:
        assert fix["max_abs_node_diff"] == 0.0 and fix["max_abs_weight_diff"] <= 4e-18


def _sto3g(zeta):
    base = [(0.444635, 0.109818), (0.535328, 0.405771), (0.154329, 2.22766)]
    prims = [(c, e * zeta ** 2) for c, e in base]
    cs = B.norm_coeff("S", [p[0] for p in prims], [p[1] for p in prims])
    return B.CGF(tuple(zip(cs, [p[1] for p in prims])), "S")


def test_h2_sto3g_textbook_integrals_and_energy():
    atoms = [B.AtomData((0.0, 0.0, 0.0), [_sto3g(1.24)], 1.0, "H"),
             B.AtomData((0.0, 0.0, 1.4), [_sto3g(1.24)], 1.0, "H")]
    fb = B.flatten(atoms)
    ob = O.OracleBasis(fb)
    s, t, eri = ob.overlap(False), ob.kinetic(), ob.eri_canonical(False)
    assert s[1] == pytest.approx(0.6593, abs=1e-4)
    assert t[0] == pytest.approx(0.7600, abs=1e-4) and t[1] == pytest.approx(0.2365, abs=1e-4)
    # (11|11), (11|12), (11|22), (12|12)
    np.testing.assert_allclose([eri[0], eri[1], eri[2], eri[3]], [0.7746, 0.4441, 0.5697, 0.2970], atol=1e-4)
    r = O.scf(fb, O.SCFOptions.baseline(direct=False))
    assert r.energy == pytest.approx(-1.1167, abs=1e-4)


def test_heh_cation_sto3g_textbook_energy():
    atoms = [B.AtomData((0.0, 0.0, 0.0), [_sto3g(2.0925)], 2.0, "He"),
             B.AtomData((0.0, 0.0, 1.4632), [_sto3g(1.24)], 1.0, "H")]
    r = O.scf(B.flatten(atoms), O.SCFOptions.reference())
    assert r.energy == pytest.approx(-2.860662, abs=2e-6)
