"""The oracle with d shells (6-31G*): direct and stored-ERI Fock builds agree,
the d components keep the reference's per-component normalisation, and the
SCF energies of the two screening paths match."""
import numpy as np

import oracle as O
from gbhf import basis as B, molecules as M


def test_d_shell_components_and_normalisation():
    fb = B.flatten(M.water_atoms("6-31g*", "text"))
    assert fb.n_cgf == 19
    lx = [tuple(int(v) for v in r) for r in fb.cgf_lxyz[9:15]]
    assert lx == [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]
    # normCoeff: Dxx carries 1/sqrt(3) of Dxy's primitive normalisation
    off = np.concatenate([[0], np.cumsum(fb.cgf_nprim)])
    c = [fb.prim_coef[off[i]] for i in range(9, 15)]
    assert abs(c[1] / c[0] - np.sqrt(3.0)) < 1e-13 and abs(c[3] / c[0] - 1.0) < 1e-13


def test_d_direct_equals_stored_fock():
    fb = B.flatten(M.water_atoms("6-31g*", "text"))
    ob = O.OracleBasis(fb)
    rng = np.random.default_rng(5)
    d = rng.standard_normal((fb.n_cgf, fb.n_cgf)) * 0.2
    d = O.square_to_tri(d + d.T)
    h = ob.hcore(False)
    f_direct, _ = ob.fock_direct(h, d, 0.0)
    np.testing.assert_allclose(f_direct, O.fock_canonical(h, d, ob.eri_canonical(False)), rtol=0, atol=1e-12)


def test_d_scf_energy():
    fb = B.flatten(M.water_atoms("6-31g*", "text"))
    e = O.scf(fb, O.SCFOptions.baseline()).energy
    assert abs(e - (-76.0104960432639)) < 1e-9
    assert abs(O.scf(fb, O.SCFOptions.baseline(guess="sad")).energy - e) < 1e-9
