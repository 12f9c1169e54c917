"""Flat layouts and index maps (NumericalTools/LinearAlgebra.hs:240-316,
HartreeFock/HartreeFock.hs:153-181) and the oracle's internal consistency."""
import numpy as np
import pytest

import oracle as O
from conftest import golden
from gbhf import basis as B, molecules as M


def canonical_keys(n):
    """calcIntegrals' enumeration (HartreeFock.hs:171-181), literally."""
    out = []
    for i in range(n):
        for j in range(i, n):
            for k in range(i, n):
                for l in range(k, n):
                    if O.sort_keys([i, j, k, l]) == [i, j, k, l]:
                        out.append((i, j, k, l))
    return out


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 9])
def test_canonical_order_and_index(n):
    keys = canonical_keys(n)
    p = n * (n + 1) // 2
    assert len(keys) == p * (p + 1) // 2
    for pos, k in enumerate(keys):
        assert O.canonical_index(n, *k) == pos
        assert O.four_index_to_flat(n, list(k)) == pos


@pytest.mark.parametrize("n", [1, 2, 5, 8])
def test_flat_index_roundtrip(n):
    idx = 0
    for i in range(n):
        for j in range(i, n):
            assert O.index_dim2_to_flat(n, i, j) == idx == O.index_dim2_to_flat(n, j, i)
            assert O.index_flat_to_dim2(n, idx) == (i, j)
            idx += 1
    assert O.dim_triang(idx) == n


def test_sort_keys_symmetry():
    rng = np.random.default_rng(0)
    for _ in range(200):
        k = list(rng.integers(0, 6, size=4))
        s = O.sort_keys(k)
        i, j, kk, l = k
        for perm in ([j, i, kk, l], [i, j, l, kk], [kk, l, i, j], [l, kk, j, i]):
            assert O.sort_keys(perm) == s


def test_water_fixture_regression():
    g = golden("water_sto3g.json")
    for variant in ("shipped", "text"):
        fb = B.flatten(M.water_atoms("sto-3g", variant))
        ob = O.OracleBasis(fb)
        for ref, key in ((True, "reference"), (False, "exact")):
            np.testing.assert_allclose(ob.overlap(ref), g[variant][key]["overlap"], rtol=0, atol=1e-14)
            np.testing.assert_allclose(ob.hcore(ref), g[variant][key]["hcore"], rtol=0, atol=1e-13)
            np.testing.assert_allclose(ob.eri_canonical(ref), g[variant][key]["eri"], rtol=0, atol=1e-14)
        assert O.scf(fb, O.SCFOptions.reference()).energy == pytest.approx(
            g[variant]["energy_reference_driver"], abs=1e-10)


def test_reference_quirks_present():
    """S_ii = 1.0 only in the reference preset; the shipped SP exponents are 1.0."""
    fb = B.flatten(M.water_atoms("sto-3g", "shipped"))
    assert np.all(fb.prim_exp[3:12] == 1.0)
    ob = O.OracleBasis(B.flatten(M.water_atoms("sto-3g", "text")))
    s_ref, s_ex = ob.overlap(True), ob.overlap(False)
    diag = [O.index_dim2_to_flat(7, i, i) for i in range(7)]
    assert np.all(s_ref[diag] == 1.0)
    assert not np.all(s_ex[diag] == 1.0)
    assert np.max(np.abs(s_ex[diag] - 1.0)) < 1e-4


def test_direct_fock_matches_stored_eri_fock():
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g", index=7))   # (H2O)2, 26 functions
    ob = O.OracleBasis(fb)
    n = fb.n_cgf
    rng = np.random.default_rng(3)
    d = rng.standard_normal((n, n)) * 0.1
    d = O.square_to_tri(d + d.T)
    h = ob.hcore(False)
    f_stored = O.fock_canonical(h, d, ob.eri_canonical(False))
    f_direct, stats = ob.fock_direct(h, d, 0.0)
    np.testing.assert_allclose(f_direct, f_stored, rtol=0, atol=1e-12)
    f_screened, st2 = ob.fock_direct(h, d, 1e-12)
    np.testing.assert_allclose(f_screened, f_stored, rtol=0, atol=1e-9)
    assert st2[2] >= 0 and st2[0] <= stats[0]


def test_cluster_energies_fixture():
    g = golden("clusters.json")
    for name, rec in g.items():
        if "batch_index" not in rec:
            continue   # (H2O)16 takes minutes on the CPU; the GPU tests check it
        fb = B.flatten(M.cluster_atoms("batch256", rec["basis"], index=rec["batch_index"]))
        r = O.scf(fb, O.SCFOptions.baseline())
        assert r.energy == pytest.approx(rec["energy"], abs=1e-9)


def test_shell_grouping():
    ob = O.OracleBasis(B.flatten(M.water_atoms("6-31g", "text")))
    sh = ob.shells()
    # O: s6, s3, p3, s1, p1 ; H: s3, s1 (x2)
    assert list(sh["L"]) == [0, 0, 1, 0, 1, 0, 0, 0, 0]
    assert list(sh["nprim"]) == [6, 3, 3, 1, 1, 3, 1, 3, 1]
    assert list(sh["ncomp"]) == [1, 1, 3, 1, 3, 1, 1, 1, 1]
